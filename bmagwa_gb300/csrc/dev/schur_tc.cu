// The exact per-SNP conditional marginal likelihood (Schur complement scan).
//
// For every chain's current model (columns X, prior precisions, upper Cholesky
// factor U of X'X + diag(inv), v = U^-T X'y, S = nu s2 + y'y - v'v) and every
// single term x = x_t(j) of every SNP outside the model, the change of the
// model's log marginal likelihood from adding x with the chain's shared prior
// precision inv_t:
//
//   u = U^-T X'x,  d2 = x'x + inv_t - u'u,  w = (x'y - u'v) / sqrt(d2)
//   dLML = 1/2 log inv_t - 1/2 log d2 - (n + nu)/2 (log(S - w^2) - log S)
//
// which is Model::update_likelihood_on_add (src/model.hpp:432-506) applied to
// each candidate without changing the model.  X'x is exact: the genotype
// columns' part is a tcgen05 GEMM of the 0/1/2 codings (products <= 4, sums
// below 2^24 for n below 4,194,304, exact in FP32), the covariate part comes
// from the exact genotype counts and fixed-point sums.  The triangular solve
// and the rest are FP64.
#include <algorithm>
#include <cstdio>

#include "tc_mainloop.cuh"

namespace {

constexpr int SC_EPI = 8;                    // epilogue warps
constexpr int SC_THREADS = 192 + 32 * SC_EPI;
constexpr int SC_KMAX = 128;                 // model columns (covariates + terms) supported

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v)
{
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

// dLML of adding term `term` of SNP j to chain c's current model; g holds X'x
// in the model's column order and is overwritten with u = U^-T X'x
__device__ double schur_unit(const DevConst& K, int c, uint64_t j, int term, double* g)
{
  const DevModel& M = K.cur[c];
  const int k = M.xcols;
  const double* U = M.l;
  for (int i = 0; i < k; ++i) {
    const double* col = U + (size_t)i * (i + 1) / 2;
    double s = g[i];
    for (int r = 0; r < i; ++r) s -= col[r] * g[r];
    g[i] = s / col[i];
  }
  double uu = 0, uv = 0;
  for (int i = 0; i < k; ++i) {
    uu += g[i] * g[i];
    uv += g[i] * M.v[i];
  }
  const DevPheno& P = K.ph[K.pheno_of[c]];
  const double inv_t = K.ch[c].inv_t2a2[term];
  const double xxc = (double)term_cross_same(P.cnt, j, term, term);
  const size_t nv = K.m_e > 1 ? K.m_e : 1;
  const int64_t* gs = P.gsum + (size_t)j * nv * 2;
  const double xy = (double)((long long)coefH(term) * gs[0] + (long long)coefR(term) * gs[1]) * ldexp(1.0, -P.sy);
  const double d2 = xxc + inv_t - uu;
  if (!(d2 > 0)) return -INFINITY;
  const double lcc = sqrt(d2);
  const double w = (xy - uv) / lcc;
  const double S = M.syx;
  return 0.5 * log(inv_t) - log(lcc) + P.minus_n_plus_nu_2 * (log(S - w * w) - log(S));
}

}  // namespace

// B rows: chain c's model genotype column r (r < its term count) at row
// c KB + r as bf16 0/1/2 codings over n_pad individuals, zero rows after it.
extern "C" __global__ void __launch_bounds__(256)
bmg_schur_cols_kernel(DevConst K, uint32_t KB, uint16_t* bm)
{
  const uint32_t row = blockIdx.x, c = row / KB, r = row % KB;
  const DevModel& M = K.cur[c];
  const int me = K.m_e;
  const int kg = M.xcols - me;
  uint16_t* dst = bm + (size_t)row * K.n_pad;
  if ((int)r >= kg) {
    for (uint64_t i = threadIdx.x; i < K.n_pad; i += blockDim.x) dst[i] = 0;
    return;
  }
  const uint32_t snp = M.xc_snp[me + r];
  const int term = M.xc_type[me + r];
  const uint8_t* codes = K.geno + (size_t)snp * K.gs;
  for (uint64_t i = threadIdx.x; i < K.n_pad; i += blockDim.x) {
    const int v = (i < K.n) ? term_value((codes[i >> 2] >> ((i & 3) * 2)) & 3, term) : 0;
    dst[i] = v == 0 ? 0 : (v == 1 ? 0x3F80 : 0x4000);
  }
}

extern "C" __global__ void __launch_bounds__(SC_THREADS, 1)
bmg_schur_tc_kernel(DevConst K, TcParams P, uint32_t KB, uint32_t n_terms, double* out,
                    const __grid_constant__ CUtensorMap map_b, const __grid_constant__ CUtensorMap map_g)
{
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  __shared__ TcCtl ctl;
  __shared__ int epi_ok;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const uint32_t ct = P.chains_tile;
  const uint32_t my_tiles = (P.tiles > blockIdx.x) ? (P.tiles - blockIdx.x + gridDim.x - 1) / gridDim.x : 0;
  const uint32_t tmem = tc_setup(P, ctl, SC_EPI);

  if (warp < 6) {
    tc_main_roles(P, ctl, smem, tmem, my_tiles, map_b, map_g);
  } else {
    // warp w reads TMEM lanes 32 (w % 4) .. +31 = rows of the tile; the two
    // warps of a quarter split the tile's chains
    const uint32_t e = warp - 6;
    const uint32_t quarter = warp & 3, part = e >> 2, nparts = SC_EPI / 4;
    const uint32_t row = quarter * 32 + lane;
    const uint32_t sl = row / P.tpad, q = row % P.tpad;
    const int term = P.term_of_row[q];
    const uint32_t c_lo = part * ct / nparts, c_hi = (part + 1) * ct / nparts;
    const int me = K.m_e;
    double g[SC_KMAX];
    for (uint32_t i = 0; i < my_tiles; ++i) {
      const uint32_t tile = blockIdx.x + i * gridDim.x;
      const uint32_t snp0 = (tile % P.m_tiles) * P.snps_per_tile;
      const uint32_t chain0 = (tile / P.m_tiles) * ct;
      const uint32_t b = i % P.n_acc, u = i / P.n_acc;
      if (e == 0) {
        bool ok = false;
        if (lane == 0) ok = !ctl.abort_flag && mbar_wait(&ctl.acc_full[b], u & 1, P.wait_limit);
        ok = __shfl_sync(0xffffffffu, ok, 0);
        if (lane == 0) {
          epi_ok = ok;
          if (!ok) ctl.abort_flag = 1;
        }
      }
      named_bar_sync(1, 32 * SC_EPI);
      if (!epi_ok) break;
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint64_t j = (uint64_t)snp0 + sl;
      const bool live_row = term >= 0 && j < K.p;
      for (uint32_t cl = c_lo; cl < c_hi; ++cl) {
        const uint32_t c = chain0 + cl;
        if (c >= K.n_chains) break;  // uniform across the warp
        const int kg = K.cur[c].xcols - me;
        __syncwarp();  // the TMEM loads are warp-wide; rows that skipped rejoin here
        // the chain's X'x entries of the genotype columns: exact integers
        for (int ch = 0; ch < kg; ch += 16) {
          float v[16];
          tmem_ld16(tmem + ((quarter * 32) << 16) + b * TC_ACC_COLS + cl * KB + ch, v);
#pragma unroll
          for (int t = 0; t < 16; ++t)
            if (ch + t < kg) g[me + ch + t] = (double)__float2int_rn(v[t]);
        }
        if (!live_row) continue;
        double& o = out[((size_t)c * K.p + j) * n_terms + q];
        if ((K.inbits[(size_t)c * ((K.p + 31) / 32) + (j >> 5)] >> (j & 31)) & 1u) {
          o = NAN;
          continue;
        }
        // covariate entries: the constant from the counts, the others from
        // the fixed-point sums
        const DevPheno& P = K.ph[K.pheno_of[c]];
        g[0] = (double)term_sum(P.cnt, j, term);
        for (int r = 1; r < me; ++r) {
          const int64_t* gs = P.gsum + ((size_t)j * me + r) * 2;
          g[r] = (double)((long long)coefH(term) * gs[0] + (long long)coefR(term) * gs[1]) * ldexp(1.0, -K.se[r]);
        }
        o = schur_unit(K, (int)c, j, term, g);
      }
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      __syncwarp();
      if (lane == 0) mbar_arrive(&ctl.acc_empty[b]);
    }
  }
  if (tc_teardown(ctl, tmem) && tid == 0) atomicExch(&K.ch[0].error, BMG_DERR_TIMEOUT);
}

// ----------------------------------------------------------------- host side

// Plan and launch.  Returns 0, or a step number on failure; 100 when a model
// is wider than the kernel supports.
extern "C" int bmg_schur_launch(const DevConst* K, const int* xcols, uint16_t** bm, size_t* bm_cap, double* out,
                                cudaStream_t stream)
{
  const uint32_t C = K->n_chains, me = K->m_e;
  uint32_t kg_max = 1;
  for (uint32_t c = 0; c < C; ++c) {
    if (xcols[c] > SC_KMAX) return 100;
    kg_max = std::max<uint32_t>(kg_max, (uint32_t)std::max(0, xcols[c] - (int)me));
  }
  const uint32_t KB = ((kg_max + 15) / 16) * 16;
  if (KB > TC_ACC_COLS || K->n >= (1u << 22) || K->n_pad % TC_BK != 0) return 1;
  TcParams P;
  const uint32_t T = K->n_terms;
  P.tpad = T <= 1 ? 1 : (T <= 2 ? 2 : 4);
  P.snps_per_tile = TC_BM / P.tpad;
  for (uint32_t u = 0; u < 4; ++u) P.term_of_row[u] = (u < T) ? K->term_of[u] : -1;
  P.k_chunks = K->n_pad / TC_BK;
  P.a_bytes = 2 * TC_A_SUB_BYTES;  // A in shared memory: the accumulators may take all 512 columns
  P.a_tmem = 0;
  P.a_stages = 0;
  P.n_acc = 2;
  P.acc_cols = TC_ACC_COLS;
  P.pk_bytes = P.snps_per_tile * (TC_BK / 4);
  P.chains_tile = std::max(1u, std::min(C, TC_ACC_COLS / KB));
  P.n_mma = P.chains_tile * KB;
  P.b_bytes = P.n_mma * TC_BK * 2;  // two 128-byte-swizzled boxes of 64 individuals
  P.stage_bytes = ((P.b_bytes + P.a_bytes + P.pk_bytes + 1023) / 1024) * 1024;
  P.xr_bytes = 0;
  P.b_rows_per_tile = P.chains_tile * KB;
  P.stages = 0;
  for (uint32_t st = TC_MAX_STAGES; st >= 2 && !P.stages; --st)
    if ((size_t)st * P.stage_bytes + 1024 <= 227 * 1024 - 9 * 1024) P.stages = st;
  if (!P.stages) return 2;
  tc_set_rings(P, P.stages);
  P.m_tiles = (uint32_t)((K->p + P.snps_per_tile - 1) / P.snps_per_tile);
  P.n_tiles = (C + P.chains_tile - 1) / P.chains_tile;
  P.tiles = P.m_tiles * P.n_tiles;
  // B: the model columns of every chain
  const size_t need = (size_t)C * KB * K->n_pad;
  if (*bm_cap < need) {
    if (*bm) cudaFree(*bm);
    *bm = nullptr;
    *bm_cap = 0;
    if (cudaMalloc(bm, need * sizeof(uint16_t)) != cudaSuccess) return 3;
    *bm_cap = need;
  }
  bmg_schur_cols_kernel<<<C * KB, 256, 0, stream>>>(*K, KB, *bm);
  if (cudaGetLastError() != cudaSuccess) return 4;
  auto enc = encode_fn();
  if (!enc) return 5;
  CUtensorMap mb, mg;
  {
    cuuint64_t dims[2] = {K->n_pad, (cuuint64_t)C * KB};
    cuuint64_t strides[1] = {(cuuint64_t)K->n_pad * 2};
    cuuint32_t box[2] = {TC_BK_SUB, P.n_mma};
    cuuint32_t es[2] = {1, 1};
    if (enc(&mb, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, (void*)*bm, dims, strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
            CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
      return 6;
  }
  {
    cuuint64_t dims[2] = {K->gs, K->p};
    cuuint64_t strides[1] = {K->gs};
    cuuint32_t box[2] = {TC_BK / 4, P.snps_per_tile};
    cuuint32_t es[2] = {1, 1};
    if (enc(&mg, CU_TENSOR_MAP_DATA_TYPE_UINT8, 2, (void*)K->geno, dims, strides, box, es,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
      return 7;
  }
  const size_t smem = (size_t)P.stages * P.stage_bytes + 1024;
  static size_t configured = 0;
  if (configured < smem) {
    if (cudaFuncSetAttribute(bmg_schur_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
        cudaSuccess)
      return 8;
    configured = smem;
  }
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (sms <= 0) sms = 1;
  const unsigned grid = (unsigned)std::min<uint32_t>(P.tiles, (uint32_t)sms);
  bmg_schur_tc_kernel<<<grid, SC_THREADS, smem, stream>>>(*K, P, KB, T, out, mb, mg);
  return cudaGetLastError() == cudaSuccess ? 0 : 9;
}
