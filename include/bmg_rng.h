/*
 * bmg_rng.h -- the random stream shared by the GPU sampler and the CPU oracle.
 *
 * The reference draws every random number of a chain from one sequential
 * generator (src/rand.hpp:174-186: boost::mt19937 feeding uniform_01,
 * normal_distribution and gamma_distribution).  Its Boost version is not
 * pinned, so the bit stream of a historical bmagwa binary cannot be
 * reproduced.  This header defines the stream instead, identically for host
 * C/C++ and CUDA device code, so that the GPU chain and the CPU oracle consume
 * the same numbers in the same order:
 *
 *   - engine: Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random
 *     numbers: as easy as 1, 2, 3", SC'11), keyed by (chain seed, 0x424d4741).
 *   - every logical draw (one uniform, one normal, one gamma variate) takes the
 *     next 64-bit "slot" of the chain; a draw that needs several raw words uses
 *     sub-counters of its own slot.  Draw k of a chain is therefore a pure
 *     function of (seed, k), which lets a p-wide scan draw per-SNP variates in
 *     parallel at known slots.
 *   - uniform_01: 53-bit double in [0, 1).
 *   - normal: Box-Muller (Box & Muller 1958), cosine branch only.
 *   - gamma(shape a): Marsaglia & Tsang (2000), "A simple method for generating
 *     gamma variables", ACM TOMS 26(3); for a < 1 the boost U^(1/a) of the same
 *     paper.  Attempts are bounded (BMG_GAMMA_MAX_TRIES); a stream that runs
 *     out returns NaN so device code can flag it instead of spinning.
 */
#ifndef BMG_RNG_H_
#define BMG_RNG_H_

#include <stdint.h>
#include <math.h>

#if defined(__CUDACC__)
#define BMG_RNG_FN __host__ __device__ __forceinline__
#else
#define BMG_RNG_FN static inline
#endif

#define BMG_RNG_KEY1 0x424d4741u        /* second key word of every chain */
#define BMG_RNG_TAG 0x6d676221u         /* fourth counter word of every block */
#define BMG_GAMMA_MAX_TRIES 64u
#define BMG_GAMMA_BOOST_SUB 0x80000000u /* sub-counter of the a<1 boost uniform */

typedef struct bmg_rng {
  uint32_t key0;  /* chain seed */
  uint32_t key1;
  uint64_t slot;  /* index of the next logical draw */
} bmg_rng_t;

BMG_RNG_FN void bmg_rng_init(bmg_rng_t* r, uint32_t seed)
{
  r->key0 = seed;
  r->key1 = BMG_RNG_KEY1;
  r->slot = 0;
}

BMG_RNG_FN void bmg_mulhilo32(uint32_t a, uint32_t b, uint32_t* hi, uint32_t* lo)
{
  uint64_t p = (uint64_t)a * (uint64_t)b;
  *hi = (uint32_t)(p >> 32);
  *lo = (uint32_t)p;
}

/* Philox4x32-10 of a 128-bit counter under a 64-bit key: ten rounds of two
   32x32->64 multiplications, the key bumped by the Weyl constants between
   rounds (the published algorithm; its known-answer vectors are checked on
   the CPU). */
BMG_RNG_FN void bmg_philox4x32_10(const uint32_t ctr[4], uint32_t key0, uint32_t key1, uint32_t out[4])
{
  uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
  uint32_t k0 = key0, k1 = key1;
  for (int round = 0; round < 10; ++round) {
    uint32_t hi0, lo0, hi1, lo1;
    bmg_mulhilo32(0xD2511F53u, c0, &hi0, &lo0);
    bmg_mulhilo32(0xCD9E8D57u, c2, &hi1, &lo1);
    uint32_t n0 = hi1 ^ c1 ^ k0;
    uint32_t n2 = hi0 ^ c3 ^ k1;
    c0 = n0; c1 = lo1; c2 = n2; c3 = lo0;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

/* One block of a chain's stream: counter (slot, sub, tag). */
BMG_RNG_FN void bmg_rng_block(uint32_t key0, uint32_t key1, uint64_t slot,
                              uint32_t sub, uint32_t out[4])
{
  const uint32_t ctr[4] = {(uint32_t)slot, (uint32_t)(slot >> 32), sub, BMG_RNG_TAG};
  bmg_philox4x32_10(ctr, key0, key1, out);
}

/* 53 random bits from two words, scaled into [0, 1). */
BMG_RNG_FN double bmg_u53(uint32_t a, uint32_t b)
{
  uint64_t m = ((uint64_t)(a >> 5) << 26) | (uint64_t)(b >> 6);
  return (double)m * (1.0 / 9007199254740992.0);
}

/* 32 random bits scaled into the open interval (0, 1). */
BMG_RNG_FN double bmg_u32open(uint32_t a)
{
  return ((double)a + 0.5) * (1.0 / 4294967296.0);
}

BMG_RNG_FN double bmg_uniform01_at(uint32_t key0, uint32_t key1, uint64_t slot)
{
  uint32_t w[4];
  bmg_rng_block(key0, key1, slot, 0u, w);
  return bmg_u53(w[0], w[1]);
}

BMG_RNG_FN double bmg_uniform01(bmg_rng_t* r)
{
  return bmg_uniform01_at(r->key0, r->key1, r->slot++);
}

/* Box-Muller on one block: u1 in (0,1], u2 in [0,1). */
BMG_RNG_FN double bmg_box_muller(uint32_t w0, uint32_t w1, uint32_t w2, uint32_t w3)
{
  double u1 = 1.0 - bmg_u53(w0, w1);
  double u2 = bmg_u53(w2, w3);
  return sqrt(-2.0 * log(u1)) * cos(6.283185307179586476925286766559 * u2);
}

BMG_RNG_FN double bmg_normal_at(uint32_t key0, uint32_t key1, uint64_t slot)
{
  uint32_t w[4];
  bmg_rng_block(key0, key1, slot, 0u, w);
  return bmg_box_muller(w[0], w[1], w[2], w[3]);
}

BMG_RNG_FN double bmg_normal(bmg_rng_t* r)
{
  return bmg_normal_at(r->key0, r->key1, r->slot++);
}

/* Gamma(shape a, scale 1) drawn from the sub-counters of one slot. */
BMG_RNG_FN double bmg_gamma_at(uint32_t key0, uint32_t key1, uint64_t slot, double a)
{
  double boost = 1.0;
  double shape = a;
  if (!(a > 0.0)) return NAN;
  if (a < 1.0) {
    uint32_t w[4];
    bmg_rng_block(key0, key1, slot, BMG_GAMMA_BOOST_SUB, w);
    boost = pow(bmg_u53(w[0], w[1]) , 1.0 / a);
    shape = a + 1.0;
  }
  double d = shape - 1.0 / 3.0;
  double c = 1.0 / sqrt(9.0 * d);
  for (uint32_t sub = 0; sub < BMG_GAMMA_MAX_TRIES; ++sub) {
    uint32_t w[4];
    bmg_rng_block(key0, key1, slot, sub, w);
    /* the normal comes from words 0,1 (radius) and word 2 (angle) */
    double u1 = 1.0 - bmg_u53(w[0], w[1]);
    double u2 = bmg_u32open(w[2]);
    double x = sqrt(-2.0 * log(u1)) * cos(6.283185307179586476925286766559 * u2);
    double v = 1.0 + c * x;
    if (v <= 0.0) continue;
    v = v * v * v;
    double u = bmg_u32open(w[3]);
    double x2 = x * x;
    if (u < 1.0 - 0.0331 * x2 * x2) return d * v * boost;
    if (log(u) < 0.5 * x2 + d * (1.0 - v + log(v))) return d * v * boost;
  }
  return NAN;
}

BMG_RNG_FN double bmg_gamma(bmg_rng_t* r, double a)
{
  return bmg_gamma_at(r->key0, r->key1, r->slot++, a);
}

#endif /* BMG_RNG_H_ */
