// CPU check of the scan's register decode (bmagwa_gb300/csrc/dev/decode_bf16.h):
// every code byte under every term coding against the codings written out
// directly.  Prints the number of mismatching 16-bit values.
#include <cstdint>
#include <cstdio>

#include "../bmagwa_gb300/csrc/dev/decode_bf16.h"

// the coding of a 2-bit code under term t (0 A, 1 H, 2 D, 3 R; -1 none)
static int coding(int code, int term)
{
  if (term < 0) return 0;
  const int g = code == 2 ? 1 : (code == 3 ? 2 : 0);
  switch (term) {
    case 0: return g;
    case 1: return g == 1;
    case 2: return g > 0;
    default: return g == 2;
  }
}

static uint32_t bf16_of(int v) { return v == 0 ? 0 : (v == 1 ? 0x3F80 : 0x4000); }

int main()
{
  long bad = 0;
  for (int term = -1; term < 4; ++term) {
    int value[4];
    for (int c = 0; c < 4; ++c) value[c] = term < 0 ? -1 : coding(c, term);
    const DecTab t = dec_tab(value);
    for (uint32_t b = 0; b < 256; ++b) {
      uint32_t o0, o1;
      dec_byte(b, t, o0, o1);
      const uint32_t got[4] = {o0 & 0xFFFF, o0 >> 16, o1 & 0xFFFF, o1 >> 16};
      for (int i = 0; i < 4; ++i)
        if (got[i] != bf16_of(coding((b >> (2 * i)) & 3, term))) ++bad;
    }
  }
  std::printf("mismatches %ld\n", bad);
  return bad != 0;
}
