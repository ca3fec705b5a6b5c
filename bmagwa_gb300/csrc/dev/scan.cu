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
    if (need) rb_epilogue(K, c, j, acc);
  }
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

// Rebuild the dd_add prefix of every chain whose proposal weights changed.
extern "C" __global__ void __launch_bounds__(1024)
bmg_rebuild_kernel(DevConst K, int force)
{
  __shared__ long long part[1024];
  const int c = blockIdx.x;
  if (!force && !K.ch[c].rebuild) return;
  rebuild_chain(K, c, part, K.ch + c);
}
