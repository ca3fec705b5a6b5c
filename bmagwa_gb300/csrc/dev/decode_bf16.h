// Packed 2-bit genotype codes -> bf16 codings with register arithmetic only
// (no tables in memory), for the A operand of the tensor-core scans.
//
// One byte of PLINK codes holds four individuals (code c_i in bits 2i, 2i+1).
// Spread: t = (b | b << 12) & 0x000F000F puts c0 c1 in bits 0-3 and c2 c3 in
// bits 16-19; (t | t << 6) & 0x03030303 leaves c_i alone in byte i.  Then
// s = t * 0x11 + 0x04040404 makes byte i the two selector nibbles
// (c_i + 4, c_i), so a byte permute of the 8-byte table {ty : tx} with
// selector s (low 16 bits) yields [lo(c0), hi(c0), lo(c1), hi(c1)]: the bf16
// codings of individuals 0 and 1 as one 32-bit word, and s >> 16 those of
// individuals 2 and 3.  tx holds the high byte of the coding of each code,
// ty the low byte (bf16 0, 1, 2 = 0x0000, 0x3F80, 0x4000).
//
// The header compiles as CUDA device code and as plain C++ (the CPU check
// compares it with the codings of every byte and term).
#ifndef BMG_DECODE_BF16_H_
#define BMG_DECODE_BF16_H_

#include <stdint.h>

#ifdef __CUDACC__
#define DEC_FN __host__ __device__ __forceinline__
#else
#define DEC_FN inline
#endif

// byte n of the result = byte ((s >> 4n) & 7) of the 8 bytes {y : x}
DEC_FN uint32_t dec_byte_perm(uint32_t x, uint32_t y, uint32_t s)
{
#if defined(__CUDA_ARCH__)
  return __byte_perm(x, y, s);
#else
  const uint64_t v = ((uint64_t)y << 32) | x;
  uint32_t r = 0;
  for (int n = 0; n < 4; ++n) r |= (uint32_t)((v >> (8 * ((s >> (4 * n)) & 7))) & 0xFF) << (8 * n);
  return r;
#endif
}

// the tables of a term from its coding of the four codes (values 0, 1, 2);
// value[c] < 0 gives zeros (rows beyond a SNP's terms)
struct DecTab {
  uint32_t x, y;
};

DEC_FN DecTab dec_tab(const int* value)
{
  DecTab t = {0, 0};
  for (int c = 0; c < 4; ++c) {
    const int v = value[c];
    const uint32_t hi = v == 1 ? 0x3F : (v == 2 ? 0x40 : 0);
    const uint32_t lo = v == 1 ? 0x80 : 0;
    t.x |= hi << (8 * c);
    t.y |= lo << (8 * c);
  }
  return t;
}

// the bf16 codings of the four individuals of code byte b: o0 = individuals
// 0, 1; o1 = individuals 2, 3 (first individual in the low half)
DEC_FN void dec_byte(uint32_t b, DecTab t, uint32_t& o0, uint32_t& o1)
{
  uint32_t s = (b | (b << 12)) & 0x000F000Fu;
  s = (s | (s << 6)) & 0x03030303u;
  s = s * 0x11u + 0x04040404u;
  o0 = dec_byte_perm(t.x, t.y, s);
  o1 = dec_byte_perm(t.x, t.y, s >> 16);
}

#endif
