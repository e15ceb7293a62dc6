// Host-side accuracy check of the double-float arithmetic of the mixed path
// (nhqg_gb300/csrc/df64.cuh), run by tests/test_df64_host.py.  The same
// operator code runs here with plain IEEE FP32 operations (compiled without
// FP contraction) as on the device with the _rn intrinsics; results are
// compared with long-double references.  Prints the worst errors and exits
// non-zero if a bound is exceeded.
#include <cmath>
#include <cstdio>
#include <random>

#include "df64.cuh"

using nhqg::dfl;

static long double ld(dfl a) { return (long double)a.hi + (long double)a.lo; }

int main() {
  std::mt19937_64 g(11);
  std::uniform_real_distribution<double> u(-1.0, 1.0);
  auto rnd = [&](int span) { return u(g) * std::ldexp(1.0, (int)(u(g) * span)); };
  // bounds: a sum within 2^-46 of |a| + |b|; a product or fma within 2^-44 of
  // |a b| (+ |c|) -- pairs straight from the truncating FP64 split carry a low
  // word up to one unit of the high word's last place, so the three FP32
  // roundings of the product's error term reach 3 x 2^-46
  const double two46 = std::ldexp(1.0, -46), two44 = std::ldexp(1.0, -44);
  double w_add = 0, w_mul = 0, w_fma = 0, w_in = 0, w_round = 0;
  long bad = 0;
  for (int i = 0; i < 2000000; ++i) {
    const double xa = rnd(40), xb = (i % 3 == 0) ? -xa * (1.0 + 1e-9 * u(g)) : rnd(40), xc = rnd(40);
    const dfl a = nhqg::df_from_double(xa), b = nhqg::df_from_double(xb), c = nhqg::df_from_double(xc);
    // FP64 -> double-float split and back
    const double ein = std::fabs((double)(ld(a) - (long double)xa)) / std::fabs(xa);
    w_in = std::fmax(w_in, ein / two46);
    const double back = nhqg::df_to_double(a);
    w_round = std::fmax(w_round, std::fabs(back - xa) / std::fabs(xa) / two46);
    // sum: error bounded relative to |a| + |b| (cancellation included)
    const long double s_ex = ld(a) + ld(b);
    const double e_add = std::fabs((double)(ld(a + b) - s_ex)) / (double)(std::fabs(ld(a)) + std::fabs(ld(b)));
    w_add = std::fmax(w_add, e_add / two46);
    // product: relative error
    const long double p_ex = ld(a) * ld(b);
    w_mul = std::fmax(w_mul, std::fabs((double)((ld(a * b) - p_ex) / p_ex)) / two44);
    // fused multiply-add: relative to |a b| + |c|
    const long double f_ex = ld(a) * ld(b) + ld(c);
    const double e_fma = std::fabs((double)(ld(nhqg::fma(a, b, c)) - f_ex)) /
                         (double)(std::fabs(p_ex) + std::fabs(ld(c)));
    w_fma = std::fmax(w_fma, e_fma / two44);
  }
  // float -> double widening is exact for normal floats, 0 below 2^-126
  for (int i = 0; i < 200000; ++i) {
    const float f = (float)rnd(120);
    const double want = (std::fabs(f) < std::ldexp(1.0f, -126)) ? 0.0 : (double)f;
    if (nhqg::f2d_bits(f) != want) ++bad;
  }
  std::printf("worst errors in units of the bound: split %.3f, round trip %.3f, add %.3f, mul %.3f, fma %.3f; "
              "widening mismatches %ld\n", w_in, w_round, w_add, w_mul, w_fma, bad);
  return (w_in <= 1.0 && w_round <= 1.0 && w_add <= 1.0 && w_mul <= 1.0 && w_fma <= 1.0 && bad == 0) ? 0 : 1;
}
