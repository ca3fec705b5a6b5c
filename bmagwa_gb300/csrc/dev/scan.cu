// The p-wide Rao-Blackwellised scan (src/sampler.cpp:32-261 and the proposal
// update :739-810) and the dd_add prefix rebuild.
//
// Products x_j' r are exact: r is a fixed-point integer vector and genotype
// codings are small integers, so both scan implementations (SIMT here, the
// tensor-core GEMM in scan_tc.cu) produce identical int64 sums.  The
// epilogue turns them into the reference's single-SNP Bayes factors.
#include <math.h>

#include "rb_epilogue.cuh"

// SIMT scan: a warp per (SNP, batch of 32 chains); lane = chain.
// The residual is read as int64 in individual-major order resid_t[i * C + c].
extern "C" __global__ void __launch_bounds__(256)
bmg_scan_simt_kernel(DevConst K, const int64_t* resid_t)
{
  const int lane = threadIdx.x & 31;
  const uint64_t warps = (uint64_t)gridDim.x * (blockDim.x >> 5);
  const uint64_t wid = (uint64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const uint32_t C = K.n_chains;
  const uint32_t nb = (C + 31) / 32;
  for (uint64_t task = wid; task < K.p * nb; task += warps) {
    uint64_t j = task / nb;
    int c = (int)(task % nb) * 32 + lane;
    bool live = c < (int)C;
    bool need = live && (K.rb[live ? c : 0].do_scan != 0);
    long long acc[4] = {0, 0, 0, 0};
    const uint8_t* row = K.geno + j * (size_t)K.gs;
    if (__any_sync(FULL_MASK, need)) {
      for (uint64_t i = 0; i < K.n; ++i) {
        int code = (row[i >> 2] >> ((i & 3) * 2)) & 3;
        if (code == 0) continue;
        long long R = live ? resid_t[i * C + c] : 0;
        int g = (code == 2) ? 1 : 2;
        acc[0] += g * R;                 // A
        if (g == 1) acc[1] += R;         // H
        acc[2] += R;                     // D
        if (g == 2) acc[3] += R;         // R
      }
    }
    if (need) {
      if (rb_fast_ok(K) && rb_plain(K, c, j)) {
        double lo;
        const double pr = rb_fast_pr(K, c, j, acc[K.types[0]], &lo);
        rb_store1(K, c, j, pr, lo);
      } else {
        rb_epilogue(K, c, j, acc);
      }
    }
  }
}

// out[i] = the scan's table-driven exp of a[i], |a[i]| <= 700 (self-test).
extern "C" __global__ void bmg_exp_selftest_kernel(const double* a, double* out, uint64_t n)
{
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
    out[i] = bmg_exp_tab(a[i]);
}

// Transpose the move kernel's residuals (chains x n_pad) to individual-major.
extern "C" __global__ void bmg_resid_transpose_kernel(DevConst K, int64_t* resid_t)
{
  uint64_t total = K.n * (uint64_t)K.n_chains;
  for (uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; t < total;
       t += (uint64_t)gridDim.x * blockDim.x) {
    uint64_t i = t / K.n_chains, c = t % K.n_chains;
    resid_t[t] = K.resid[c * K.n_pad + i];
  }
}

// Rebuild the dd_add prefix of every chain whose proposal weights changed
// (or of all chains with force), in two passes over tiles of
// BMG_REBUILD_TILE in-order positions: tile sums, then each tile's exclusive
// prefix written with its offset.  The weights and their order are those of
// rebuild_chain (common.cuh).
extern "C" __global__ void __launch_bounds__(256)
bmg_rebuild_sums_kernel(DevConst K, int force)
{
  __shared__ long long red[8];
  const uint32_t t = blockIdx.x, c = blockIdx.y;
  const bool active = force || K.ch[c].rebuild;
  if (t == 0 && threadIdx.x == 0) K.rebuild_active[c] = active;
  if (!active) return;
  const uint64_t p = K.p, q0 = (uint64_t)t * BMG_REBUILD_TILE;
  const uint64_t q1 = min(p, q0 + BMG_REBUILD_TILE);
  const double* pp = K.p_prop + (size_t)c * p;
  const uint32_t* ib = K.inbits + (size_t)c * ((p + 31) / 32);
  const double sc = ldexp(1.0, K.qs);
  long long sum = 0;
  for (uint64_t q = q0 + threadIdx.x; q < q1; q += blockDim.x) {
    const uint32_t snp = (uint32_t)K.inv[q];
    if (!((ib[snp >> 5] >> (snp & 31)) & 1u)) sum += __double2ll_rn(fmax(pp[q], K.q_add_min) * sc);
  }
  sum = warp_sum_ll(sum);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = sum;
  __syncthreads();
  if (threadIdx.x == 0) {
    long long tot = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) tot += red[w];
    K.tile_sums[(size_t)c * gridDim.x + t] = tot;
  }
}

extern "C" __global__ void __launch_bounds__(256)
bmg_rebuild_write_kernel(DevConst K)
{
  constexpr int PER = BMG_REBUILD_TILE / 256;  // consecutive positions per thread
  __shared__ long long part[256];
  __shared__ long long base_sh;
  const uint32_t t = blockIdx.x, c = blockIdx.y, tiles = gridDim.x;
  if (!K.rebuild_active[c]) return;
  const int tid = threadIdx.x;
  const uint64_t p = K.p;
  // offset of this tile: the sum of the earlier tiles' sums
  if (tid < 32) {
    long long o = 0;
    for (uint32_t u = tid; u < t; u += 32) o += K.tile_sums[(size_t)c * tiles + u];
    o = warp_sum_ll(o);
    if (tid == 0) base_sh = o;
  }
  const double* pp = K.p_prop + (size_t)c * p;
  const uint32_t* ib = K.inbits + (size_t)c * ((p + 31) / 32);
  const double sc = ldexp(1.0, K.qs);
  const uint64_t q0 = (uint64_t)t * BMG_REBUILD_TILE + (uint64_t)tid * PER;
  long long w[PER];
  long long mine = 0;
#pragma unroll
  for (int r = 0; r < PER; ++r) {
    const uint64_t q = q0 + r;
    long long v = 0;
    if (q < p) {
      const uint32_t snp = (uint32_t)K.inv[q];
      if (!((ib[snp >> 5] >> (snp & 31)) & 1u)) v = __double2ll_rn(fmax(pp[q], K.q_add_min) * sc);
    }
    w[r] = v;
    mine += v;
  }
  part[tid] = mine;
  __syncthreads();
  for (int o = 1; o < 256; o <<= 1) {
    long long v = (tid >= o) ? part[tid - o] : 0;
    __syncthreads();
    part[tid] += v;
    __syncthreads();
  }
  long long run = base_sh + part[tid] - mine;
  int64_t* cadd = K.cadd + (size_t)c * (p + 1);
#pragma unroll
  for (int r = 0; r < PER; ++r) {
    const uint64_t q = q0 + r;
    if (q < p) cadd[q] = run;
    run += w[r];
  }
  // the zero state of the new base: this tile's share of the bitmap words
  const uint64_t nwords = (p + 31) / 32;
  uint32_t* bb = K.basebits + (size_t)c * nwords;
  for (uint64_t wd = (uint64_t)t * (BMG_REBUILD_TILE / 32) + tid; wd < min(nwords, (uint64_t)(t + 1) * (BMG_REBUILD_TILE / 32));
       wd += blockDim.x)
    bb[wd] = ib[wd];
  if (t == tiles - 1 && tid == 255) {
    cadd[p] = run;
    K.ch[c].cadd_total = run;
    K.ch[c].n_pend = 0;
    K.ch[c].rebuild = 0;
  }
}
