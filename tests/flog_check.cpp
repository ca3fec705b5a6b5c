// CPU check of the move kernel's table-driven logarithm (bmagwa_gb300/csrc/
// dev/flog.h) against long double: prints the largest error in ulps of the
// result over seeded random arguments across the double range, near 1 and
// at the table's break points.  Built with -ffp-contract=off by
// tests/test_df64.py (the FMAs are explicit).
#include <cfloat>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <random>

#define __device__
#define __forceinline__ inline
using std::fma;
using std::log;
#include "../bmagwa_gb300/csrc/dev/flog.h"

static double ulps(double got, double x)
{
  const long double ref = logl((long double)x);
  const double r = (double)ref;
  const double u = r == 0 ? DBL_MIN : std::nextafter(std::fabs(r), INFINITY) - std::fabs(r);
  return (double)(fabsl((long double)got - ref) / u);
}

int main()
{
  std::mt19937_64 g(777);
  std::uniform_real_distribution<double> ue(-1000, 1000), u01(0, 1), near(-1e-3, 1e-3);
  double worst = 0, worst_x = 0, worst_near1 = 0;
  for (int i = 0; i < 2000000; ++i) {
    const double x = std::exp2(ue(g)) * (1 + u01(g));
    const double e = ulps(flog(x), x);
    if (e > worst) { worst = e; worst_x = x; }
  }
  for (int i = 0; i < 1000000; ++i) {
    const double x = 1 + near(g);
    const double e = ulps(flog(x), x);
    if (e > worst_near1) worst_near1 = e;
  }
  double worst_unit = 0;
  std::uniform_real_distribution<double> u0515(0.5, 2.0);
  for (int i = 0; i < 2000000; ++i) {
    const double x = u0515(g);
    const double e = ulps(flog(x), x);
    if (e > worst_unit) worst_unit = e;
  }
  double worst_break = 0;
  for (int j = 0; j < 256; ++j)
    for (int k = -3; k <= 3; ++k) {
      const double x = std::nextafter(1.0 + j / 256.0, k < 0 ? 0.0 : 2.0);
      for (int s = -2; s <= 2; ++s) {
        const double xs = std::ldexp(x, s * 7);
        const double e = ulps(flog(xs), xs);
        if (e > worst_break) worst_break = e;
      }
    }
  const bool special = flog(0.0) == -INFINITY && std::isnan(flog(-1.0)) && flog(INFINITY) == INFINITY &&
                       flog(1.0) == 0.0 && std::fabs(flog(4.9e-324) - std::log(4.9e-324)) == 0;
  std::printf("random %.3f\nnear1 %.3f\nunit %.3f\nbreaks %.3f\nspecial %d\n", worst, worst_near1, worst_unit,
              worst_break, special ? 1 : 0);
  std::fprintf(stderr, "worst at %a\n", worst_x);
  return 0;
}
