// The pair scans' CCD yes/no (ccd_hits, ccd2d.hpp) against the full test (ccd_happens, the
// reference's ballBallCCDCollisionHappens with its square root and divisions): the same answer on
// disc pairs like a pile's, on quadratics built with roots at a hair's breadth from 0 and 1, on
// random bit patterns (NaN, infinities, subnormals, huge values) and on a grid of special values.
// Compiled with -ffp-contract=off, as the device code is with -fmad=false.  Exit status 0 = pass.
#include "ccd2d.hpp"

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <random>

int main(int argc, char** argv) {
  const long n_cases = argc > 1 ? std::atol(argv[1]) : 2000000;
  std::mt19937_64 g(20260412);
  std::uniform_real_distribution<double> u(-1.0, 1.0);
  long bad = 0, n = 0;
  auto check = [&](double c0, double c1, double c2) {
    const bool a = sg::ccd_happens(c0, c1, c2, nullptr), b = sg::ccd_hits(c0, c1, c2);
    ++n;
    if (a != b) {
      if (bad < 10) std::printf("mismatch c0=%a c1=%a c2=%a: ccd_happens %d ccd_hits %d\n", c0, c1, c2, a, b);
      ++bad;
    }
  };
  for (long k = 0; k < n_cases; ++k) {
    const double ra = 0.04 + 0.01 * (u(g) + 1.0), rb = 0.04 + 0.01 * (u(g) + 1.0);
    const double dx = u(g) * 0.15, dy = u(g) * 0.15;
    const double s = (k % 3 == 0) ? 1e-3 : (k % 3 == 1 ? 1e-6 : 1e-1);
    const double ex = u(g) * s, ey = u(g) * s, rs = ra + rb;
    check((dx * dx + dy * dy) - rs * rs, 2.0 * (dx * ex + dy * ey), ex * ex + ey * ey);
  }
  for (long k = 0; k < n_cases; ++k) {
    const double c2 = std::ldexp(1.0 + 0.5 * u(g), (int)(u(g) * 60));
    double r0 = 1.0 + u(g) * std::ldexp(1.0, -(int)(10 + 45 * (0.5 + 0.5 * u(g))));
    double r1 = r0 + std::fabs(u(g)) * std::ldexp(1.0, -(int)(50 * (0.5 + 0.5 * u(g))));
    if (k & 1) {
      const double t = -r1;
      r1 = -r0;
      r0 = t;
    }
    const double c1 = -c2 * (r0 + r1), c0 = c2 * r0 * r1;
    check(c0, c1, c2);
    check(c0, -c1, c2);
    check(c0, std::nextafter(c1, 0.0), c2);
  }
  for (long k = 0; k < n_cases; ++k) {
    std::uint64_t b[3] = {g(), g(), g()};
    double c[3];
    std::memcpy(c, b, sizeof c);
    check(c[0], c[1], std::fabs(c[2]));
    check(std::fabs(c[0]), c[1], std::fabs(c[2]));
  }
  const double sp[] = {0.0, -0.0, 1e-320, -1e-320, 0x1p-500, 0x1p500, 0x1.fffffffffffffp499, 0x1p-501, 0x1p501,
                       1.0, -1.0, 2.0, 0.5, -0.5, 1e300, -1e300, INFINITY, -INFINITY, NAN};
  for (double a : sp)
    for (double b : sp)
      for (double c : sp) check(a, b, std::fabs(c));
  std::printf("%ld cases, %ld mismatches\n", n, bad);
  return bad == 0 ? 0 : 1;
}
