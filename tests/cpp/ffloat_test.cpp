// The float-float pairs of the FP64-precision disc sweeps (ffloat.hpp) on the host: the split of a
// double keeps 48 bits, hi + lo is exact in FP64, and sums, products and a long accumulation stay
// within small multiples of 2^-48 of their operands' magnitudes, against long double arithmetic.
// Compiled with -ffp-contract=off, as the device code is built without contraction.
// Exit status 0 = pass.
#include "ffloat.hpp"

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <random>

using sg::FF;

static long g_bad = 0;

static void expect(bool ok, const char* what, double a, double b, long double err, long double bound) {
  if (!ok) {
    if (g_bad < 10)
      std::printf("%s: a=%.17g b=%.17g err=%Lg bound=%Lg\n", what, a, b, err, bound);
    ++g_bad;
  }
}

int main(int argc, char** argv) {
  const long n = argc > 1 ? std::atol(argv[1]) : 1000000;
  std::mt19937_64 g(7);
  std::uniform_real_distribution<double> u(-1.0, 1.0);
  std::uniform_int_distribution<int> ex(-30, 30);
  const long double e48 = std::ldexp(1.0L, -48), e44 = std::ldexp(1.0L, -44);
  for (long k = 0; k < n; ++k) {
    const double a = std::ldexp(u(g), ex(g)), b = (k % 4 == 0) ? -a * (1.0 + std::ldexp(u(g), -30))
                                                                : std::ldexp(u(g), ex(g));
    const FF fa = sg::ff_split(a), fb = sg::ff_split(b);
    const double va = sg::ff_value(fa), vb = sg::ff_value(fb);
    // split: 48 bits, and hi + lo exact in FP64
    expect(std::fabs((long double)va - a) <= e48 * std::fabs(a), "split", a, 0, std::fabs((long double)va - a),
           e48 * std::fabs(a));
    expect((long double)fa.hi + (long double)fa.lo == (long double)va, "value exact", a, 0, 0, 0);
    const long double m = std::fmax(std::fabs(va), std::fabs(vb));
    // sum and difference
    const long double s = (long double)va + (long double)vb;
    const long double es = std::fabs((long double)sg::ff_value(sg::ff_add(fa, fb)) - s);
    expect(es <= e44 * m, "add", a, b, es, e44 * m);
    const long double d = (long double)va - (long double)vb;
    const long double ed = std::fabs((long double)sg::ff_value(sg::ff_sub(fa, fb)) - d);
    expect(ed <= e44 * m, "sub", a, b, ed, e44 * m);
    // product
    const long double p = (long double)va * (long double)vb;
    const long double ep = std::fabs((long double)sg::ff_value(sg::ff_mul(fa, fb)) - p);
    expect(ep <= e44 * std::fabs(p), "mul", a, b, ep, e44 * std::fabs(p));
    // pair + float
    const float f = (float)b;
    const long double sf = (long double)va + (long double)f;
    const long double ef = std::fabs((long double)sg::ff_value(sg::ff_add_f(fa, f)) - sf);
    expect(ef <= e44 * std::fmax(std::fabs(va), std::fabs((double)f)), "add_f", a, f, ef,
           e44 * std::fmax(std::fabs(va), std::fabs((double)f)));
  }
  // A velocity accumulated over many impulse increments, as in a long solve: v += m * p.
  for (int trial = 0; trial < 20; ++trial) {
    FF v = sg::ff_split(u(g) * 0.05);
    long double vl = sg::ff_value(v);
    const FF mi = sg::ff_split(800.0 * (0.5 + 0.5 * std::fabs(u(g))));
    const long double ml = sg::ff_value(mi);
    long double vmax = std::fabs(vl);
    const int steps = 20000;
    for (int k = 0; k < steps; ++k) {
      const FF p = sg::ff_split(u(g) * 1e-6);
      v = sg::ff_add(v, sg::ff_mul(mi, p));
      vl += ml * (long double)sg::ff_value(p);
      vmax = std::fmax(vmax, std::fabs(vl));
    }
    const long double err = std::fabs((long double)sg::ff_value(v) - vl);
    expect(err <= steps * e44 * vmax, "accumulation", 0, 0, err, steps * e44 * vmax);
  }
  std::printf("%ld checks failed\n", g_bad);
  return g_bad == 0 ? 0 : 1;
}
