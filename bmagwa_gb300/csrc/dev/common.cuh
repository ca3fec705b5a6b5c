// Device helpers shared by the libbmg kernels.
#ifndef BMG_DEV_COMMON_CUH_
#define BMG_DEV_COMMON_CUH_

#include <stdint.h>
#include <cuda_runtime.h>

#include "state.h"

#define FULL_MASK 0xffffffffu

__device__ __forceinline__ int lane_id() { return threadIdx.x & 31; }
__device__ __forceinline__ int warp_id() { return threadIdx.x >> 5; }

__device__ __forceinline__ double warp_sum_d(double v)
{
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(FULL_MASK, v, o);
  return v;
}

__device__ __forceinline__ long long warp_sum_ll(long long v)
{
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(FULL_MASK, v, o);
  return v;
}

__device__ __forceinline__ int warp_sum_i(int v)
{
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(FULL_MASK, v, o);
  return v;
}

__device__ __forceinline__ double shfl_d(double v, int src)
{
  return __shfl_sync(FULL_MASK, v, src);
}

// 2-bit PLINK code of individual i in a genotype row
__device__ __forceinline__ int geno_code(const uint8_t* row, uint64_t i)
{
  return (row[i >> 2] >> ((i & 3) * 2)) & 3;
}

// a genotype 0/1/2 in term coding t (A, H, D, R; src/genotype_tables.hpp)
__device__ __forceinline__ int gval_term(int g, int t)
{
  return t == 0 ? g : (t == 1 ? (g == 1) : (t == 2 ? (g > 0) : (g == 2)));
}

// imputed genotype of a missing call from the cumulative counts of the SNP's
// calls (DataModel::sample_missing, src/data_model.cpp:78-103, one uniform
// through Utils::sample_discrete_naive, src/utils.cpp:46-57)
__device__ __forceinline__ int miss_draw(const double* mp, double u)
{
  const double r = u * mp[2];
  return r < mp[0] ? 0 : (r < mp[1] ? 1 : 2);
}

// genotype value of a term coding from a 2-bit code (00->0, 10->1, 11->2;
// src/data.cpp:36 and src/genotype_tables.hpp).  Missing codes never reach
// the device path (they are rejected at load).
__device__ __forceinline__ int term_value(int code, int term)
{
  int g = (code == 2) ? 1 : (code == 3 ? 2 : 0);
  switch (term) {
    case 0: return g;
    case 1: return g == 1;
    case 2: return g > 0;
    default: return g == 2;
  }
}

// Coefficients of the H = [g==1] and R = [g==2] indicator planes in a term
// coding: A = H + 2R, H = H, D = H + R, R = R.
__device__ __forceinline__ int coefH(int term) { return term == 3 ? 0 : 1; }
__device__ __forceinline__ int coefR(int term) { return term == 0 ? 2 : (term == 1 ? 0 : 1); }

// sum over individuals of a term's values from the genotype counts
__device__ __forceinline__ int64_t term_sum(const int32_t* cnt, uint64_t snp, int term)
{
  int64_t n1 = cnt[2 * snp], n2 = cnt[2 * snp + 1];
  return coefH(term) * n1 + coefR(term) * n2;
}

// cross product of two codings of the same SNP: sum_i x_t(g_i) x_u(g_i)
__device__ __forceinline__ int64_t term_cross_same(const int32_t* cnt, uint64_t snp, int t, int u)
{
  int64_t n1 = cnt[2 * snp], n2 = cnt[2 * snp + 1];
  return (int64_t)coefH(t) * coefH(u) * n1 + (int64_t)coefR(t) * coefR(u) * n2;
}

__device__ __forceinline__ uint64_t ld_u64(const uint8_t* p) { return *(const uint64_t*)p; }


// Rebuild the dd_add prefix of chain c with the calling CTA (all threads):
// weights in the in-order position order of the reference's proposal tree
// (src/discrete_distribution.hpp:217-314), zero for SNPs in the current
// model, exclusive prefix sums in fixed point (weight * 2^qs).  The totals
// go to `chain` (the chain's state in global or shared memory).
__device__ inline void rebuild_chain(const DevConst& K, int c, long long* part, DevChain* chain)
{
  const int tid = threadIdx.x, nth = blockDim.x;
  const uint64_t p = K.p;
  const uint64_t per = (p + nth - 1) / nth;
  const uint64_t q0 = min(p, (uint64_t)tid * per), q1 = min(p, q0 + per);
  const double* pp = K.p_prop + (size_t)c * p;
  const uint32_t* ib = K.inbits + (size_t)c * ((p + 31) / 32);
  const double sc = ldexp(1.0, K.qs);
  long long sum = 0;
  for (uint64_t q = q0; q < q1; ++q) {
    uint32_t snp = (uint32_t)K.inv[q];
    bool z = (ib[snp >> 5] >> (snp & 31)) & 1u;
    if (!z) sum += __double2ll_rn(fmax(pp[q], K.q_add_min) * sc);
  }
  __syncthreads();
  part[tid] = sum;
  __syncthreads();
  for (int o = 1; o < nth; o <<= 1) {
    long long v = (tid >= o) ? part[tid - o] : 0;
    __syncthreads();
    part[tid] += v;
    __syncthreads();
  }
  long long run = part[tid] - sum;
  int64_t* cadd = K.cadd + (size_t)c * (p + 1);
  for (uint64_t q = q0; q < q1; ++q) {
    cadd[q] = run;
    uint32_t snp = (uint32_t)K.inv[q];
    bool z = (ib[snp >> 5] >> (snp & 31)) & 1u;
    if (!z) run += __double2ll_rn(fmax(pp[q], K.q_add_min) * sc);
  }
  uint32_t* bb = K.basebits + (size_t)c * ((p + 31) / 32);
  for (uint64_t w = tid; w < (p + 31) / 32; w += nth) bb[w] = ib[w];
  __syncthreads();
  if (tid == nth - 1) {
    cadd[p] = part[nth - 1];
    chain->cadd_total = part[nth - 1];
    chain->n_pend = 0;
    chain->rebuild = 0;
  }
  __syncthreads();
}

#endif
