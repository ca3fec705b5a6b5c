/* Host check of the random stream header (include/bmg_rng.h), compiled as C:
 * the Philox4x32-10 block on the published known-answer counters, then
 * moments of each variate the sampler draws, as "name value" lines. */
#include <stdio.h>

#include "bmg_rng.h"

static void kat(const char* name, uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, uint32_t k0, uint32_t k1)
{
  const uint32_t ctr[4] = {c0, c1, c2, c3};
  uint32_t out[4];
  bmg_philox4x32_10(ctr, k0, k1, out);
  printf("%s %08x%08x%08x%08x\n", name, out[0], out[1], out[2], out[3]);
}

int main(void)
{
  kat("kat_zero", 0, 0, 0, 0, 0, 0);
  kat("kat_ones", 0xffffffffu, 0xffffffffu, 0xffffffffu, 0xffffffffu, 0xffffffffu, 0xffffffffu);
  kat("kat_pi", 0x243f6a88u, 0x85a308d3u, 0x13198a2eu, 0x03707344u, 0xa4093822u, 0x299f31d0u);

  const long N = 4000000;
  bmg_rng_t r;
  bmg_rng_init(&r, 1234u);
  double s1 = 0, s2 = 0, lo = 1, hi = 0;
  for (long i = 0; i < N; ++i) {
    double u = bmg_uniform01(&r);
    s1 += u;
    s2 += u * u;
    if (u < lo) lo = u;
    if (u > hi) hi = u;
  }
  printf("uniform_mean %.10g\nuniform_var %.10g\nuniform_min %.10g\nuniform_max %.10g\n", s1 / N,
         s2 / N - (s1 / N) * (s1 / N), lo, hi);

  double m[5] = {0, 0, 0, 0, 0};
  for (long i = 0; i < N; ++i) {
    double x = bmg_normal(&r), p = 1;
    for (int k = 1; k <= 4; ++k) {
      p *= x;
      m[k] += p;
    }
  }
  printf("normal_m1 %.10g\nnormal_m2 %.10g\nnormal_m3 %.10g\nnormal_m4 %.10g\n", m[1] / N, m[2] / N, m[3] / N,
         m[4] / N);

  const double shapes[6] = {0.3, 0.5, 1.0, 2.5, 10.0, 100.0};
  long nan_count = 0;
  for (int k = 0; k < 6; ++k) {
    double a = shapes[k], g1 = 0, g2 = 0;
    for (long i = 0; i < N / 4; ++i) {
      double g = bmg_gamma(&r, a);
      if (g != g) {
        ++nan_count;
        continue;
      }
      g1 += g;
      g2 += g * g;
    }
    double mean = g1 / (N / 4), var = g2 / (N / 4) - mean * mean;
    printf("gamma_mean_%g %.10g\ngamma_var_%g %.10g\n", a, mean, a, var);
  }
  printf("gamma_nan %ld\n", nan_count);
  /* the slot of draw k is k: the same draw from a fresh stream at slot 7 */
  bmg_rng_t a, b;
  bmg_rng_init(&a, 99u);
  bmg_rng_init(&b, 99u);
  for (int i = 0; i < 7; ++i) bmg_normal(&a);
  b.slot = 7;
  printf("slot_addressable %d\n", bmg_gamma(&a, 2.5) == bmg_gamma(&b, 2.5));
  return 0;
}
