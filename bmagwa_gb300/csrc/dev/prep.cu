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

// Exact fixed-point sums of the phenotype (v = 0) and of covariate v (v >= 1)
// over the heterozygous and the homozygous-alternate individuals of every
// SNP: gsum[(j * nv + v) * 2 + {0, 1}].  A term's product with the vector is
// then coefH * H-sum + coefR * R-sum, exactly the sum over individuals of
// x_t(g_i) * vec_i that Model::update_add needs for X'y and X'E
// (src/model.hpp:432-506).  One warp per SNP; each lane takes whole bytes
// (4 individuals); the vectors are staged through shared memory in chunks.
#define GSUM_CHUNK 2048
extern "C" __global__ void __launch_bounds__(256)
bmg_gsum_kernel(const uint8_t* geno, uint64_t n, uint64_t p, uint32_t gs, const int64_t* yint,
                const int64_t* eint, uint32_t nv, int64_t* gsum)
{
  __shared__ int64_t vec[GSUM_CHUNK];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const uint64_t snps_per_block = blockDim.x >> 5;
  for (uint64_t base = (uint64_t)blockIdx.x * snps_per_block; base < p; base += (uint64_t)gridDim.x * snps_per_block) {
    const uint64_t j = base + warp;
    const uint8_t* row = geno + (j < p ? j : 0) * gs;
    for (uint32_t v = 0; v < nv; ++v) {
      const int64_t* src = (v == 0) ? yint : eint + (size_t)v * n;
      long long sh = 0, sr = 0;
      for (uint64_t c0 = 0; c0 < n; c0 += GSUM_CHUNK) {
        const uint64_t len = min((uint64_t)GSUM_CHUNK, n - c0);
        __syncthreads();
        for (uint64_t i = threadIdx.x; i < len; i += blockDim.x) vec[i] = src[c0 + i];
        __syncthreads();
        if (j < p) {
          for (uint64_t b = lane; b < (len + 3) / 4; b += 32) {
            uint32_t byte = row[(c0 >> 2) + b];
#pragma unroll
            for (int q = 0; q < 4; ++q) {
              const uint64_t i = 4 * b + q;
              const int code = (byte >> (2 * q)) & 3;
              if (i < len) {
                if (code == 2) sh += vec[i];
                else if (code == 3) sr += vec[i];
              }
            }
          }
        }
      }
      sh = warp_sum_ll(sh);
      sr = warp_sum_ll(sr);
      if (j < p && lane == 0) {
        gsum[(j * nv + v) * 2] = sh;
        gsum[(j * nv + v) * 2 + 1] = sr;
      }
    }
  }
}

// Several phenotypes: #het and #hom-alt of every SNP among the individuals of
// every sample (mask2: 01 in the 2-bit slot of each individual of sample k),
// cnt[(k p + j) 2 + {0, 1}].  One warp per (SNP, sample).
extern "C" __global__ void __launch_bounds__(256)
bmg_mask_counts_kernel(const uint8_t* geno, uint32_t gs, uint64_t p, const uint64_t* mask2, uint32_t n_samples,
                       int32_t* cnt)
{
  const int lane = threadIdx.x & 31;
  const uint64_t warps = (uint64_t)gridDim.x * (blockDim.x >> 5);
  const uint64_t nw64 = gs / 8;
  // SNP-major: consecutive warps take the samples of one SNP, so its row is
  // read from memory once and from cache by the others (the masks, gs / 4
  // bytes per sample, stay in L2)
  for (uint64_t q = (uint64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); q < p * n_samples; q += warps) {
    const uint64_t j = q / n_samples, k = q % n_samples, t = k * p + j;
    const uint64_t* row = reinterpret_cast<const uint64_t*>(geno + j * gs);
    const uint64_t* mk = mask2 + k * nw64;
    unsigned h = 0, r = 0;
    for (uint64_t w = lane; w < nw64; w += 32) {
      const uint64_t x = row[w], m = mk[w];
      const uint64_t hi = (x >> 1) & m, lo = x & m;
      h += __popcll(hi & ~lo);
      r += __popcll(hi & lo);
    }
    h = (unsigned)warp_sum_i((int)h);
    r = (unsigned)warp_sum_i((int)r);
    if (lane == 0) {
      cnt[t * 2] = (int32_t)h;
      cnt[t * 2 + 1] = (int32_t)r;
    }
  }
}

// The precomputed sums of every SNP within every sample from its counts
// (src/precomputed_snp_covariances.hpp:95-131; the same expressions as the
// single-sample host pass), pre[(k p + j) offset + .].
extern "C" __global__ void bmg_pre_kernel(const int32_t* cnt, uint64_t p, uint32_t n_samples, const double* n_of,
                                          int allow_mask, int ah, int offset, double* pre)
{
  for (uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; t < p * n_samples;
       t += (uint64_t)gridDim.x * blockDim.x) {
    const double n = n_of[t / p];
    const double n1 = cnt[2 * t], n2 = cnt[2 * t + 1];
    double* loc = pre + t * (uint64_t)offset;
    for (int u = 0; u < 4; ++u) {
      if (!((allow_mask >> u) & 1)) continue;
      const double ch = (u == 3) ? 0 : 1, cr = (u == 0) ? 2 : (u == 1 ? 0 : 1);
      const double xs = ch * n1 + cr * n2;
      const double xx = ch * ch * n1 + cr * cr * n2;
      *loc++ = xs;
      *loc++ = xx - xs * xs / n;
    }
    if (ah) {
      const double as = n1 + 2 * n2, hs = n1;
      *loc = n1 - as * hs / n;
    }
  }
}

// Per SNP the two precomputed sums of the scan's one-type posterior as FP32:
// out[j] = {sum x (an integer below 2^24), pre1 hi, pre1 lo, 0} with pre1 the
// centred second moment, split into a float pair (about 48 bits).
extern "C" __global__ void bmg_pre_df_kernel(const double* pre, uint64_t p, uint32_t offset, uint32_t off,
                                             float4* out)
{
  for (uint64_t j = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; j < p; j += (uint64_t)gridDim.x * blockDim.x) {
    const double* loc = pre + j * offset + off;
    const float h = (float)loc[1];
    out[j] = make_float4((float)loc[0], h, (float)(loc[1] - (double)h), 0.0f);
  }
}

// Clear the codes past the last individual in byte `last` of every row (the
// .bed format pads a row to whole bytes with unspecified bits).
extern "C" __global__ void bmg_tail_kernel(uint8_t* g, uint64_t p, uint64_t gs, uint64_t last, uint8_t keep)
{
  for (uint64_t j = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; j < p; j += (uint64_t)gridDim.x * blockDim.x)
    g[j * gs + last] &= keep;
}
