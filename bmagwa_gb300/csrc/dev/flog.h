// Natural logarithm in few FP64 instructions, for the move kernel's scalar
// path.
//
// On GB300 an FP64 instruction occupies an SM sub-partition's FP64 pipe for
// about 64 cycles whatever the number of active lanes, and the library log()
// costs about a microsecond.  flog() is a table-driven logarithm after
// Tang ("Table-driven implementation of the logarithm function in IEEE
// floating-point arithmetic", ACM TOMS 16(4), 1990) in about twelve FP64
// instructions:
//
//   x = 2^e m, m in [1, 2);  j = the top 8 fraction bits of m;
//   r_j ~ 1 / (1 + j/256) (a double from the table);  u = m r_j - 1 by one
//   FMA, so |u| < 2^-8 and u carries one rounding;
//   log x = e ln 2 - log r_j + log1p(u),
//   log1p(u) = u + u^2 (-1/2 + u/3 - u^2/4 + u^3/5 - u^4/6 + u^5/7)
//   (truncation below u^8 / 8 < 2^-67, and below 2^-59 relative to log1p u).
// Arguments within 2^-8 of 1 take u = x - 1 (exact) and no table term, so that
// the result keeps its relative accuracy where log x is small.
//
// -log r_j comes from the table as hi + lo doubles and ln 2 as a 42-bit head
// (exact times any exponent) plus a tail, so the result is within a few ulp of
// log x (checked on the host against long double by tests/test_df64.py).
// Zero, negative, subnormal, infinite and NaN arguments take log().
#ifndef BMG_FLOG_H_
#define BMG_FLOG_H_

#include <stdint.h>

#include "log_table.h"

__device__ __forceinline__ double flog(double x)
{
  if (!(x >= 2.2250738585072014e-308) || !(x <= 1.7976931348623157e308)) return log(x);
  uint64_t b;
#ifdef __CUDA_ARCH__
  b = (uint64_t)__double_as_longlong(x);
#else
  __builtin_memcpy(&b, &x, 8);
#endif
  // 1 - 2^-8 < x < 1 + 2^-8, compared as bit patterns (positive doubles
  // order as integers)
  const bool near1 = b > 0x3FEFE00000000000ull && b < 0x3FF0100000000000ull;
  const int e = near1 ? 0 : (int)((b >> 52) & 0x7FF) - 1023;
  const int j = near1 ? 0 : (int)((b >> 44) & 0xFF);
  const uint64_t mb = (b & 0x000FFFFFFFFFFFFFull) | 0x3FF0000000000000ull;
  double m;
#ifdef __CUDA_ARCH__
  m = __longlong_as_double((long long)mb);
#else
  __builtin_memcpy(&m, &mb, 8);
#endif
  const double u = near1 ? x - 1.0 : fma(m, kLogR[j], -1.0);
  const double u2 = u * u;
  const double q =
      fma(fma(fma(fma(fma(1.0 / 7.0, u, -1.0 / 6.0), u, 1.0 / 5.0), u, -0.25), u, 1.0 / 3.0), u, -0.5);
  const double p = fma(u2, q, u);
  if (near1) return p;
  const double ed = (double)e;
  const double hi = fma(ed, BMG_LN2_HI, kLogT[2 * j]);
  const double lo = fma(ed, BMG_LN2_LO, kLogT[2 * j + 1]) + p;
  return hi + lo;
}

#endif
