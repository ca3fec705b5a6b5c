// CPU check of the scan's double-float arithmetic (bmagwa_gb300/csrc/dev/
// df64.h, rb_df.h) against long double: prints the largest relative error of
// each routine and of the posterior over seeded random inputs.  Built with
// -ffp-contract=off by tests/test_df64.py.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <random>

#define __device__
#include "../bmagwa_gb300/csrc/dev/exp_table.h"
#include "../bmagwa_gb300/csrc/dev/rb_df.h"

static long double ld(dfl x) { return (long double)x.h + (long double)x.l; }

static dfl to_df(long double v)
{
  const float h = (float)v;
  return {h, (float)(v - (long double)h)};
}

static long double rel(long double got, long double ref)
{
  const long double d = fabsl(got - ref);
  return ref == 0 ? d : d / fabsl(ref);
}

int main()
{
  std::mt19937_64 g(12345);
  std::uniform_real_distribution<double> u(0.0, 1.0);
  long double e_add = 0, e_mul = 0, e_div = 0, e_rsqrt = 0, e_exp = 0, e_pr = 0, e_ll = 0;
  for (int it = 0; it < 200000; ++it) {
    const long double xa = (u(g) - 0.5) * std::pow(10.0, 8 * u(g) - 4);
    const long double xb = (u(g) - 0.3) * std::pow(10.0, 8 * u(g) - 4);
    const dfl a = to_df(xa), b = to_df(xb);
    const long double A = ld(a), B = ld(b);
    if (A + B != 0) e_add = fmaxl(e_add, rel(ld(df_add(a, b)), A + B));
    e_mul = fmaxl(e_mul, rel(ld(df_mul(a, b)), A * B));
    e_div = fmaxl(e_div, rel(ld(df_div(a, b)), A / B));
    const dfl p = to_df(fabsl(xa) + 1e-3L);
    e_rsqrt = fmaxl(e_rsqrt, rel(ld(df_rsqrt(p)), 1.0L / sqrtl(ld(p))));
    const dfl x = to_df(-60.0L + 147.0L * u(g));
    e_exp = fmaxl(e_exp, rel(ld(df_exp(x, kExp2TabF)), expl(ld(x))));
    const long long v = (long long)((u(g) - 0.5) * 9.0e18);
    e_ll = fmaxl(e_ll, rel(ld(df_from_ll(v)), (long double)v));
  }
  // the posterior on inputs shaped like a scan: n individuals, additive
  // coding, residual fixed point 2^-40, the odds spanning p_r from ~1e-20 to 1
  for (int it = 0; it < 200000; ++it) {
    const double n = 1000 + 19000 * u(g);
    const double maf = 0.05 + 0.45 * u(g);
    const double sx = std::floor(2 * maf * n);
    const double var = 2 * maf * (1 - maf) * n * (0.8 + 0.4 * u(g));
    const double itv = std::pow(10.0, 3 * u(g) - 1);
    const double mr = (u(g) - 0.5) * 1e-3;
    const double sigma2 = 0.3 + u(g);
    const double cadd = -12 - 3 * u(g);
    const double scale = std::ldexp(1.0, -40);
    const double target = 0.5 * std::sqrt(var) * (20 * u(g));  // |rx s| up to ~10 sd
    const double xr = (u(g) < 0.5 ? -1 : 1) * target * std::sqrt(var) + sx * mr;
    const long long xi = (long long)std::llround(xr / scale);
    const double pr = rb_pr_df(xi, (float)scale, (float)sx, to_df(var), to_df(mr), to_df(itv),
                               to_df(0.5L / sigma2), to_df(cadd), kExp2TabF);
    // reference: the same quantities in long double
    const long double X = (long double)xi * scale, RX = X - (long double)sx * (long double)mr;
    const long double DET = (long double)var + (long double)itv;
    const long double A = RX * RX / DET / (2.0L * sigma2) + cadd;
    const long double E = expl(A) / sqrtl(DET);
    const long double PR = E / (1 + E);
    if (pr < 0) {
      if (A >= -59.9L) e_pr = 1;  // the FP64 fallback only below -60
      continue;
    }
    e_pr = fmaxl(e_pr, rel(pr, PR));
  }
  std::printf("add %.3Le\nmul %.3Le\ndiv %.3Le\nrsqrt %.3Le\nexp %.3Le\nll %.3Le\npr %.3Le\n", e_add, e_mul, e_div,
              e_rsqrt, e_exp, e_ll, e_pr);
  return 0;
}
