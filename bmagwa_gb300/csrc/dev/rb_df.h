// The single-SNP posterior of the Rao-Blackwell scan (src/sampler.cpp:89-258,
// one effect type, shared tau2, SNP outside the model) in double-float
// arithmetic.  The same function runs in the scan kernels and in the CPU
// checks of the arithmetic.
//
// With det = x'x - (sum x)^2/n + inv_tau2 (pre1 + itv), s = det^-1/2 and
// rx = x'r - (sum x) mean(r), the log posterior odds of inclusion are
//   lo = (rx s)^2 / (2 sigma2) - log(det)/2 - slq/2 + lmp
// and p_r = exp(lo) / (1 + exp(lo)).  Here exp(lo) is evaluated as
// exp(a) s with a = (rx s)^2 / (2 sigma2) + cadd, cadd = lmp - slq/2, which
// needs no logarithm.
#ifndef BMG_RB_DF_H_
#define BMG_RB_DF_H_

#include "df64.h"

// p_r from the exact product xi = x'R (fixed point, value xi * scale, scale a
// power of two), sx = sum x (an integer below 2^24), pre1, and the chain's
// mr = mean(r), itv = inv_tau2 alpha^2, i2s = 1/(2 sigma2), cadd.  Returns 1
// when the odds exceed 2^54 (a > 87, p_r rounds to 1 in FP64; also a NaN, as
// the reference maps a non-finite exp to 1) and -1 when a < -60, which the
// caller evaluates in FP64.
DF_FN double rb_pr_df(long long xi, float scale, float sx, dfl pre1, dfl mr, dfl itv, dfl i2s, dfl cadd,
                      const float* exp_tab)
{
  dfl x = df_from_ll(xi);
  x.h = df_m(x.h, scale);
  x.l = df_m(x.l, scale);
  const dfl rx = df_add(x, df_neg(df_mul_f(mr, sx)));
  const dfl s = df_rsqrt(df_add(pre1, itv));
  const dfl t = df_mul(rx, s);
  const dfl a = df_add(df_mul(df_mul(t, t), i2s), cadd);
  if (!(a.h <= 87.0f)) return 1.0;
  if (a.h < -60.0f) return -1.0;
  const dfl e = df_mul(df_exp(a, exp_tab), s);
  return df_to_double(df_div(e, df_add_f(e, 1.0f)));
}

#endif
