// Genotype preparation on the device (src/data.cpp:324-376, src/data.cpp:403-434):
// per-SNP genotype counts, the minor-allele recode, and the missing-call
// check.  One warp per SNP; rows are read as 32-bit words of 16 individuals.
#include "common.cuh"

// counts[4*j + {0,1,2,3}] = #code00, #code10 (het), #code11, #code01 (missing)
__device__ __forceinline__ void count_word(uint32_t w, uint32_t valid_mask, unsigned* c)
{
  const uint32_t m5 = 0x55555555u;
  uint32_t lo = w & m5, hi = (w >> 1) & m5;
  uint32_t v = valid_mask & m5;
  c[0] += __popc(~hi & ~lo & v);
  c[1] += __popc(hi & ~lo & v);
  c[2] += __popc(hi & lo & v);
  c[3] += __popc(~hi & lo & v);
}

__device__ __forceinline__ uint32_t valid_bits(uint64_t n, uint64_t w)
{
  uint64_t first = w * 16;
  if (first + 16 <= n) return 0xffffffffu;
  if (first >= n) return 0u;
  uint64_t k = n - first;  // individuals in this word
  return (uint32_t)((1ull << (2 * k)) - 1);
}

// Counts, recode to minor-allele count when asked (swap codes 00 and 11 when
// the allele frequency of the current coding exceeds 0.5), counts again.
// cnt gets (#het, #hom-alt) after the recode; missing gets the missing count.
extern "C" __global__ void bmg_prep_kernel(uint8_t* geno, uint64_t n, uint64_t p, uint32_t gs,
                                           int recode, int32_t* cnt, int32_t* missing)
{
  const int lane = threadIdx.x & 31;
  const uint64_t warps = (uint64_t)gridDim.x * (blockDim.x >> 5);
  const uint64_t nw = gs / 4;
  for (uint64_t j = (uint64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); j < p; j += warps) {
    uint32_t* row = (uint32_t*)(geno + j * gs);
    unsigned c[4] = {0, 0, 0, 0};
    for (uint64_t w = lane; w < nw; w += 32) count_word(row[w], valid_bits(n, w), c);
    for (int q = 0; q < 4; ++q) c[q] = warp_sum_i((int)c[q]);
    long long ngenos = (long long)n - c[3];
    long long macount = (long long)c[1] + 2ll * c[2];
    bool swap = recode && (macount > ngenos);  // macount / (2 ngenos) > 0.5
    if (swap) {
      const uint32_t m5 = 0x55555555u;
      for (uint64_t w = lane; w < nw; w += 32) {
        uint32_t x = row[w];
        uint32_t same = ~((x >> 1) ^ x) & m5 & valid_bits(n, w);  // code 00 or 11
        row[w] = x ^ (same | (same << 1));
      }
    }
    if (lane == 0) {
      cnt[2 * j] = (int32_t)c[1];
      cnt[2 * j + 1] = (int32_t)(swap ? c[0] : c[2]);
      missing[j] = (int32_t)c[3];
    }
  }
}

extern "C" __global__ void bmg_trace_reset_kernel(DevChain* ch, int n_chains)
{
  int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c < n_chains) {
    ch[c].tr_iter = 0;
    ch[c].tr_thin = 0;
    ch[c].tr_loci = 0;
    ch[c].tr_beta = 0;
    ch[c].tr_log = 0;
  }
}
