// Double-float ("double-word") arithmetic: a value is an unevaluated sum
// hi + lo of two FP32 numbers with |lo| <= ulp(hi) / 2, giving about 44 bits
// of precision at FP32 speed.  On GB300 the FP32 pipes issue 64 times as many
// operations as the FP64 pipe, so the per-SNP posterior of the scan runs in
// this arithmetic and only the running means stay in FP64.
//
// Building blocks: Knuth's TwoSum and Dekker's FastTwoSum (D. E. Knuth, The
// Art of Computer Programming vol. 2, 4.2.2; T. J. Dekker, "A floating-point
// technique for extending the available precision", Numer. Math. 18, 1971),
// the FMA-based TwoProd, and the double-word algorithms of M. Joldes,
// J.-M. Muller and V. Popescu, "Tight and rigorous error bounds for basic
// building blocks of double-word arithmetic", ACM TOMS 44(2), 2017
// (AccurateDWPlusDW, DWTimesFP3, DWTimesDW3, DWDivDW2; relative error bounds
// 3u^2 .. 15u^2 with u = 2^-24).  Every operation rounds to nearest and must
// not be contracted or reassociated: device code uses the _rn intrinsics,
// host code (the CPU checks) is compiled with -ffp-contract=off.
//
// The header compiles as CUDA device code and as plain C++.
#ifndef BMG_DF64_H_
#define BMG_DF64_H_

#include <math.h>
#include <stdint.h>

#ifdef __CUDACC__
#define DF_FN __host__ __device__ __forceinline__
#else
#define DF_FN inline
#endif

struct dfl {
  float h, l;
};

#if defined(__CUDA_ARCH__)
DF_FN float df_a(float a, float b) { return __fadd_rn(a, b); }
DF_FN float df_s(float a, float b) { return __fsub_rn(a, b); }
DF_FN float df_m(float a, float b) { return __fmul_rn(a, b); }
DF_FN float df_f(float a, float b, float c) { return __fmaf_rn(a, b, c); }
DF_FN float df_d(float a, float b) { return __fdiv_rn(a, b); }
DF_FN float df_rsqrt_approx(float a) { return rsqrtf(a); }
#else
DF_FN float df_a(float a, float b) { return a + b; }
DF_FN float df_s(float a, float b) { return a - b; }
DF_FN float df_m(float a, float b) { return a * b; }
DF_FN float df_f(float a, float b, float c) { return fmaf(a, b, c); }
DF_FN float df_d(float a, float b) { return a / b; }
DF_FN float df_rsqrt_approx(float a) { return 1.0f / sqrtf(a); }
#endif

// s + e = a + b exactly (any magnitudes)
DF_FN dfl two_sum(float a, float b)
{
  const float s = df_a(a, b);
  const float bb = df_s(s, a);
  const float e = df_a(df_s(a, df_s(s, bb)), df_s(b, bb));
  return {s, e};
}

// s + e = a + b exactly, for |a| >= |b| (or a = 0)
DF_FN dfl fast_two_sum(float a, float b)
{
  const float s = df_a(a, b);
  return {s, df_s(b, df_s(s, a))};
}

// p + e = a b exactly (no underflow)
DF_FN dfl two_prod(float a, float b)
{
  const float p = df_m(a, b);
  return {p, df_f(a, b, -p)};
}

DF_FN dfl df_from_double(double x)
{
  const float h = (float)x;
  return {h, (float)(x - (double)h)};
}

DF_FN double df_to_double(dfl x) { return (double)x.h + (double)x.l; }

// AccurateDWPlusDW
DF_FN dfl df_add(dfl x, dfl y)
{
  const dfl s = two_sum(x.h, y.h);
  const dfl t = two_sum(x.l, y.l);
  const dfl v = fast_two_sum(s.h, df_a(s.l, t.h));
  return fast_two_sum(v.h, df_a(t.l, v.l));
}

DF_FN dfl df_neg(dfl x) { return {-x.h, -x.l}; }

// DWPlusFP
DF_FN dfl df_add_f(dfl x, float y)
{
  const dfl s = two_sum(x.h, y);
  return fast_two_sum(s.h, df_a(x.l, s.l));
}

// DWTimesFP3
DF_FN dfl df_mul_f(dfl x, float y)
{
  const dfl c = two_prod(x.h, y);
  return fast_two_sum(c.h, df_f(x.l, y, c.l));
}

// DWTimesDW3
DF_FN dfl df_mul(dfl x, dfl y)
{
  const dfl c = two_prod(x.h, y.h);
  const float tl0 = df_m(x.l, y.l);
  const float tl1 = df_f(x.h, y.l, tl0);
  const float cl2 = df_f(x.l, y.h, tl1);
  return fast_two_sum(c.h, df_a(c.l, cl2));
}

// DWDivDW2
DF_FN dfl df_div(dfl x, dfl y)
{
  const float th = df_d(x.h, y.h);
  const dfl r = df_mul_f(y, th);
  const float d = df_a(df_s(x.h, r.h), df_s(x.l, r.l));
  return fast_two_sum(th, df_d(d, y.h));
}

// 1 / sqrt(x), x > 0: the FP32 estimate y (relative error below 2^-21)
// refined with e = 1 - x y^2 (from TwoProd and DWTimesDW3) by the series
// 1/sqrt(1 - e) = 1 + e/2 + 3e^2/8 + O(e^3); the truncation is below 2^-60
DF_FN dfl df_rsqrt(dfl x)
{
  const float y = df_rsqrt_approx(x.h);
  const dfl xy2 = df_mul(x, two_prod(y, y));
  const float e = df_s(df_s(1.0f, xy2.h), xy2.l);  // 1 - xy2.h is exact (Sterbenz)
  return fast_two_sum(y, df_m(df_m(y, e), df_f(e, 0.375f, 0.5f)));
}

// exp(a) for -60 <= a.h <= 87 by Tang's method (P. T. P. Tang, ACM TOMS
// 15(2), 1989) in double-float: a = k ln2/256 + r, k = 256 m + i,
// |r| <= ln2/512; exp(a) = 2^m T_i (1 + (exp(r) - 1)) with T_i = 2^(i/256) as
// a float pair (tab[2i], tab[2i + 1]).  ln2/256 = C1 + C2 + C3 with C1 of 9
// significant bits, so k C1 is exact for |k| < 2^15, and the reduction is a
// double-float sum of exact terms (C3 k in FP32).  exp(r) - 1 =
// r + r^2/2 + r^3/6 + r^4/24 (truncation below 4e-17): r^2/2 from TwoProd,
// the cubic and quartic terms in FP32.  The result stays a normal FP32 pair
// for a >= -60.
DF_FN dfl df_exp(dfl a, const float* tab)
{
  const float C1 = 0x1.63p-9f, C2 = -0x1.bd0106p-21f, C3 = 0x1.cf79acp-48f;
  const float kf = rintf(df_m(a.h, 0x1.715476p+8f));
  const int k = (int)kf;
  dfl r = df_add_f(two_sum(a.h, -df_m(kf, C1)), a.l);  // k C1 is exact
  r = df_add(r, df_neg(two_prod(kf, C2)));
  r = df_add_f(r, df_m(-kf, C3));
  // r^2 / 2 (with the cross term r.h r.l)
  dfl q = two_prod(r.h, r.h);
  q.h = df_m(q.h, 0.5f);
  q.l = df_f(r.h, r.l, df_m(q.l, 0.5f));
  const float c34 = df_f(df_m(q.h, q.h), 1.0f / 6.0f, df_m(df_m(r.h, q.h), 1.0f / 3.0f));
  const dfl em1 = df_add_f(df_add(r, q), c34);
  const int i = k & 255, m = k >> 8;
  const dfl T = {tab[2 * i], tab[2 * i + 1]};
  const dfl y = df_add(T, df_mul(T, em1));
#if defined(__CUDA_ARCH__)
  const float sc = __int_as_float((m + 127) << 23);
#else
  const float sc = ldexpf(1.0f, m);
#endif
  return {df_m(y.h, sc), df_m(y.l, sc)};
}

// int64 -> double-float (about 48 bits of the value)
DF_FN dfl df_from_ll(long long v)
{
  const float h = (float)v;
  const long long rest = v - (long long)h;
  return {h, (float)rest};
}

#endif
